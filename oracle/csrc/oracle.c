/*
 * Plain C (OpenMP) restatement of the reference's stencil arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/ as a second oracle and by bench.py
 * as the timed CPU baseline ("port").  The product library never links it.
 *
 * Arithmetic order follows the reference's numpy verification exactly, with
 * one rounding per operation (build with -ffp-contract=off, no fast-math):
 *   hdiff  stencil_benchmarks/benchmarks_collection/stencils/base.py:284-311
 *   vadv   stencil_benchmarks/benchmarks_collection/stencils/base.py:410-473
 *   triad  stencil_benchmarks/benchmarks_collection/stream/cuda_hip.j2:158-163
 *
 * Pointers address the first interior point; strides are in elements and
 * shared by all fields (as in the reference, where every field of a stencil
 * is allocated with the same shape, layout and alignment).
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* horizontal diffusion: one k-plane per work item, lap/flx/fly rows staged  */
/* in thread-local planes so every value is computed once                    */
/* ------------------------------------------------------------------------ */
#define DEFINE_HDIFF(T, SUFFIX, FOUR)                                                  \
    int oracle_hdiff_##SUFFIX(const T* inp, const T* coeff, T* out, int64_t ni,        \
                              int64_t nj, int64_t nk, int64_t si, int64_t sj,          \
                              int64_t sk) {                                             \
        if (ni <= 0 || nj <= 0 || nk <= 0) return 0;                                   \
        const int64_t li = ni + 2, lj = nj + 2; /* lap on [-1, ni] x [-1, nj] */       \
        int failed = 0;                                                                 \
        _Pragma("omp parallel") {                                                       \
            T* lap = (T*)malloc(sizeof(T) * (size_t)(li * lj));                         \
            T* flx = (T*)malloc(sizeof(T) * (size_t)((ni + 1) * nj));                   \
            T* fly = (T*)malloc(sizeof(T) * (size_t)(ni * (nj + 1)));                   \
            if (!lap || !flx || !fly) {                                                 \
                _Pragma("omp atomic write") failed = 1;                                 \
            } else {                                                                    \
                _Pragma("omp for schedule(static)")                                     \
                for (int64_t k = 0; k < nk; ++k) {                                      \
                    const T* in = inp + k * sk;                                         \
                    for (int64_t j = -1; j <= nj; ++j)                                  \
                        for (int64_t i = -1; i <= ni; ++i) {                            \
                            const T* p = in + i * si + j * sj;                          \
                            lap[(j + 1) * li + (i + 1)] =                               \
                                FOUR * p[0] - (((p[si] + p[-si]) + p[sj]) + p[-sj]);    \
                        }                                                               \
                    /* flx at i in [-1, ni-1], j in [0, nj-1] */                        \
                    for (int64_t j = 0; j < nj; ++j)                                    \
                        for (int64_t i = -1; i < ni; ++i) {                             \
                            const T* p = in + i * si + j * sj;                          \
                            T f = lap[(j + 1) * li + (i + 2)] - lap[(j + 1) * li + (i + 1)]; \
                            flx[j * (ni + 1) + (i + 1)] = (f * (p[si] - p[0]) > 0) ? (T)0 : f; \
                        }                                                               \
                    /* fly at i in [0, ni-1], j in [-1, nj-1] */                        \
                    for (int64_t j = -1; j < nj; ++j)                                   \
                        for (int64_t i = 0; i < ni; ++i) {                              \
                            const T* p = in + i * si + j * sj;                          \
                            T f = lap[(j + 2) * li + (i + 1)] - lap[(j + 1) * li + (i + 1)]; \
                            fly[(j + 1) * ni + i] = (f * (p[sj] - p[0]) > 0) ? (T)0 : f; \
                        }                                                               \
                    for (int64_t j = 0; j < nj; ++j)                                    \
                        for (int64_t i = 0; i < ni; ++i) {                              \
                            const int64_t o = i * si + j * sj + k * sk;                 \
                            T d = ((flx[j * (ni + 1) + (i + 1)] - flx[j * (ni + 1) + i]) + \
                                   fly[(j + 1) * ni + i]) - fly[j * ni + i];            \
                            out[o] = inp[o] - coeff[o] * d;                             \
                        }                                                               \
                }                                                                       \
            }                                                                           \
            free(lap);                                                                  \
            free(flx);                                                                  \
            free(fly);                                                                  \
        }                                                                               \
        return failed ? 1 : 0;                                                          \
    }

DEFINE_HDIFF(double, f64, 4.0)
DEFINE_HDIFF(float, f32, 4.0f)

/* ------------------------------------------------------------------------ */
/* vertical advection (u component: wcon read at i+1).  One j-row of columns */
/* per work item; ccol/dcol kept in row-planes [nk][ni] so the i loop        */
/* vectorises.  tensstage is read in the forward sweep; the result goes to */
/* `out` (== tensstage for the reference's in-place update).               */
/* ------------------------------------------------------------------------ */
#define DEFINE_VADV(T, SUFFIX, DTR, QUARTER, HALF, ONE)                                  \
    int oracle_vadv_##SUFFIX(const T* stage, const T* pos, const T* tens, const T* tensstage, \
                             const T* wcon, T* out, int64_t ni, int64_t nj, int64_t nk,   \
                             int64_t si, int64_t sj, int64_t sk, int64_t wshift_i,       \
                             int64_t wshift_j) {                                          \
        if (ni <= 0 || nj <= 0) return 0;                                                \
        if (nk < 2) return 2;                                                             \
        const int64_t wsh = wshift_i * si + wshift_j * sj;                                \
        int failed = 0;                                                                   \
        _Pragma("omp parallel") {                                                         \
            T* ccol = (T*)malloc(sizeof(T) * (size_t)(nk * ni));                          \
            T* dcol = (T*)malloc(sizeof(T) * (size_t)(nk * ni));                          \
            T* data = (T*)malloc(sizeof(T) * (size_t)ni);                                 \
            if (!ccol || !dcol || !data) {                                                \
                _Pragma("omp atomic write") failed = 1;                                   \
            } else {                                                                      \
                const T dtr = DTR;                                                        \
                _Pragma("omp for schedule(static)")                                       \
                for (int64_t j = 0; j < nj; ++j) {                                        \
                    const int64_t row = j * sj;                                           \
                    /* k = 0 */                                                           \
                    for (int64_t i = 0; i < ni; ++i) {                                    \
                        const int64_t o = row + i * si;                                   \
                        T gcv = QUARTER * (wcon[o + sk + wsh] + wcon[o + sk]);            \
                        T cs = gcv * HALF;                                                \
                        T c = gcv * HALF;                                                 \
                        T bcol = dtr - c;                                                 \
                        T corr = -cs * (stage[o + sk] - stage[o]);                        \
                        T d = dtr * pos[o] + tens[o] + tensstage[o] + corr;               \
                        ccol[i] = c / bcol;                                               \
                        dcol[i] = d / bcol;                                               \
                    }                                                                     \
                    for (int64_t k = 1; k < nk - 1; ++k) {                                \
                        T* cc = ccol + k * ni;                                            \
                        T* dc = dcol + k * ni;                                            \
                        const T* cp = ccol + (k - 1) * ni;                                \
                        const T* dp = dcol + (k - 1) * ni;                                \
                        for (int64_t i = 0; i < ni; ++i) {                                \
                            const int64_t o = row + i * si + k * sk;                      \
                            T gav = -QUARTER * (wcon[o + wsh] + wcon[o]);                 \
                            T gcv = QUARTER * (wcon[o + sk + wsh] + wcon[o + sk]);        \
                            T as_ = gav * HALF;                                           \
                            T cs = gcv * HALF;                                            \
                            T acol = gav * HALF;                                          \
                            T c = gcv * HALF;                                             \
                            T bcol = dtr - acol - c;                                      \
                            T corr = -as_ * (stage[o - sk] - stage[o]) -                  \
                                     cs * (stage[o + sk] - stage[o]);                     \
                            T d = dtr * pos[o] + tens[o] + tensstage[o] + corr;           \
                            T divided = ONE / (bcol - cp[i] * acol);                      \
                            cc[i] = c * divided;                                          \
                            dc[i] = (d - dp[i] * acol) * divided;                         \
                        }                                                                 \
                    }                                                                     \
                    {                                                                     \
                        const int64_t k = nk - 1;                                         \
                        const T* cp = ccol + (k - 1) * ni;                                \
                        const T* dp = dcol + (k - 1) * ni;                                \
                        T* dc = dcol + k * ni;                                            \
                        for (int64_t i = 0; i < ni; ++i) {                                \
                            const int64_t o = row + i * si + k * sk;                      \
                            T gav = -QUARTER * (wcon[o + wsh] + wcon[o]);                 \
                            T as_ = gav * HALF;                                           \
                            T acol = gav * HALF;                                          \
                            T bcol = dtr - acol;                                          \
                            T corr = -as_ * (stage[o - sk] - stage[o]);                   \
                            T d = dtr * pos[o] + tens[o] + tensstage[o] + corr;           \
                            dc[i] = (d - dp[i] * acol) / (bcol - cp[i] * acol);           \
                        }                                                                 \
                    }                                                                     \
                    for (int64_t i = 0; i < ni; ++i) {                                    \
                        const int64_t o = row + i * si + (nk - 1) * sk;                   \
                        data[i] = dcol[(nk - 1) * ni + i];                                \
                        out[o] = dtr * (data[i] - pos[o]);                                \
                    }                                                                     \
                    for (int64_t k = nk - 2; k >= 0; --k)                                 \
                        for (int64_t i = 0; i < ni; ++i) {                                \
                            const int64_t o = row + i * si + k * sk;                      \
                            data[i] = dcol[k * ni + i] - ccol[k * ni + i] * data[i];      \
                            out[o] = dtr * (data[i] - pos[o]);                            \
                        }                                                                 \
                }                                                                         \
            }                                                                             \
            free(ccol);                                                                   \
            free(dcol);                                                                   \
            free(data);                                                                   \
        }                                                                                 \
        return failed ? 1 : 0;                                                            \
    }

DEFINE_VADV(double, f64, (3.0 / 20.0), 0.25, 0.5, 1.0)
DEFINE_VADV(float, f32, ((float)(3.0 / 20.0)), 0.25f, 0.5f, 1.0f)

/* ------------------------------------------------------------------------ */
/* STREAM triad a = b + s*c, two roundings                                   */
/* ------------------------------------------------------------------------ */
void oracle_triad_f64(double* a, const double* b, const double* c, double s, int64_t n) {
    _Pragma("omp parallel for schedule(static)")
    for (int64_t i = 0; i < n; ++i) a[i] = b[i] + s * c[i];
}
