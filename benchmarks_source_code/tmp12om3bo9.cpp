


#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iostream>

#include <errno.h>
#include <omp.h>
#ifdef __AVX__
#include <immintrin.h>
#endif


using index_t = std::int64_t;
  using vec_t = double __attribute__((vector_size(8 * sizeof(double))));
  using ivec_t = index_t __attribute__((vector_size(8 * sizeof(index_t))));

  __attribute__((always_inline)) inline vec_t loadu(const double* ptr) {
#ifdef __clang__
    ptr = (double*)__builtin_assume_aligned(ptr, sizeof(double));
    vec_t v;
    for (int i = 0; i < 8; ++i)
      v[i] = ptr[i];
    return v;
#else
  using uvec_t = double __attribute__((vector_size(8 * sizeof(double)), aligned(sizeof(double))));
  return *(uvec_t*)ptr;
#endif
  }

  __attribute__((always_inline)) inline void storeu(double* ptr, vec_t v) {
#ifdef __clang__
    ptr = (double*)__builtin_assume_aligned(ptr, sizeof(double));
    for (int i = 0; i < 8; ++i)
      ptr[i] = v[i];
#else
    using uvec_t = double __attribute__((vector_size(8 * sizeof(double)), aligned(sizeof(double))));
    *(uvec_t*)ptr = v;
#endif
  }
    __attribute__((always_inline)) inline vec_t load(const double* ptr) { return loadu(ptr); }
    __attribute__((always_inline)) inline void store(double* ptr, vec_t v) { storeu(ptr, v); }
    __attribute__((always_inline)) inline void storent(double* ptr, vec_t v) { storeu(ptr, v); }

#ifdef __clang__
  __attribute__((always_inline)) inline vec_t select(ivec_t condition, vec_t v1, vec_t v2) {
    vec_t v;
    for (int i = 0; i < 8; ++i)
      v[i] = condition[i] ? v1[i] : v2[i];
    return v;
  }
#else
  #define select(condition, v1, v2) ((condition) ? (v1) : (v2))
#endif

#ifdef __clang__
  #define shuffle(v1, v2, ...) __builtin_shufflevector(v1, v2, __VA_ARGS__)
#else
  #define shuffle(v1, v2, ...) __builtin_shuffle(v1, v2, (ivec_t){__VA_ARGS__})
#endif



#if defined(__amd64__) || defined(__x86_64__)
#include <xmmintrin.h>
#endif

static constexpr double dtr_stage = 3.0 / 20.0;
static constexpr double beta_v = 0;
static constexpr double bet_m = 0.5 * (1.0 - beta_v);
static constexpr double bet_p = 0.5 * (1.0 + beta_v);

#ifndef __clang__
#pragma omp declare simd linear(i) uniform(j, ishift, jshift, ccol, dcol, wcon, ustage, upos, utens, utensstage)
#endif
__attribute__((always_inline)) inline void forward_sweep(int i,
    const int j,
    const int ishift,
    const int jshift,
    double *__restrict__ ccol,
    double *__restrict__ dcol,
    const double *__restrict__ wcon,
    const double *__restrict__ ustage,
    const double *__restrict__ upos,
    const double *__restrict__ utens,
    const double *__restrict__ utensstage) {

    double ccol0, ccol1;
    double dcol0, dcol1;
    double ustage0, ustage1, ustage2;
    double wcon0, wcon1;
    double wcon_shift0, wcon_shift1;

    int index = i * 1 + j * 514;
    // k minimum
    {
        wcon_shift0 = wcon[index + ishift * 1 + jshift * 514 + 264196];
        wcon0 = wcon[index + 264196];
        double gcv = double(0.25) * (wcon_shift0 + wcon0);
        double cs = gcv * bet_m;

        ccol0 = gcv * bet_p;
        double bcol = dtr_stage - ccol0;

        ustage0 = ustage[index + 264196];
        ustage1 = ustage[index];
        double correction_term = -cs * (ustage0 - ustage1);
        dcol0 = dtr_stage * upos[index] + utens[index] + utensstage[index] + correction_term;

        double divided = double(1.0) / bcol;
        ccol0 = ccol0 * divided;
        dcol0 = dcol0 * divided;

        ccol[0] = ccol0;
        dcol[0] = dcol0;

        index += 264196;
    }

    // k body
    for (int k = 1; k < 80 - 1; ++k) {
        

        ccol1 = ccol0;
        dcol1 = dcol0;
        ustage2 = ustage1;
        ustage1 = ustage0;
        wcon1 = wcon0;
        wcon_shift1 = wcon_shift0;

        double gav = double(-0.25) * (wcon_shift1 + wcon1);
        wcon_shift0 = wcon[index + ishift * 1 + jshift * 514 + 264196];
        wcon0 = wcon[index + 264196];
        double gcv = double(0.25) * (wcon_shift0 + wcon0);

        double as = gav * bet_m;
        double cs = gcv * bet_m;

        double acol = gav * bet_p;
        ccol0 = gcv * bet_p;
        double bcol = dtr_stage - acol - ccol0;

        ustage0 = ustage[index + 264196];
        double correction_term = -as * (ustage2 - ustage1) - cs * (ustage0 - ustage1);
        dcol0 = dtr_stage * upos[index] + utens[index] + utensstage[index] + correction_term;

        double divided = double(1.0) / (bcol - ccol1 * acol);
        ccol0 = ccol0 * divided;
        dcol0 = (dcol0 - dcol1 * acol) * divided;

        ccol[k] = ccol0;
        dcol[k] = dcol0;

        index += 264196;
    }

    // k maximum
    {
        ccol1 = ccol0;
        dcol1 = dcol0;
        ustage2 = ustage1;
        ustage1 = ustage0;
        wcon1 = wcon0;
        wcon_shift1 = wcon_shift0;

        double gav = double(-0.25) * (wcon_shift1 + wcon1);

        double as = gav * bet_m;

        double acol = gav * bet_p;
        double bcol = dtr_stage - acol;

        double correction_term = -as * (ustage2 - ustage1);
        dcol0 = dtr_stage * upos[index] + utens[index] + utensstage[index] + correction_term;

        double divided = double(1.0) / (bcol - ccol1 * acol);
        dcol0 = (dcol0 - dcol1 * acol) * divided;

        dcol[79] = dcol0;
        ccol[79] = ccol0;
    }
}

#ifndef __clang__
#pragma omp declare simd linear(i) uniform(j, ccol, dcol, upos, utensstage)
#endif
__attribute__((always_inline)) inline void backward_sweep(int i,
    const int j,
    const double *__restrict__ ccol,
    const double *__restrict__ dcol,
    const double *__restrict__ upos,
    double *__restrict__ utensstage) {
    constexpr double dtr_stage = 3.0 / 20.0;

    double datacol;

    int index = i * 1 + j * 514 + (80 - 1) * 264196;
    // k
    {
        datacol = dcol[79];
        utensstage[index] = dtr_stage * (datacol - upos[index]);

        index -= 264196;
    }

    // k body
    for (int k = 80 - 2; k >= 0; --k) {
        datacol = dcol[k] - ccol[k] * datacol;
        utensstage[index] = dtr_stage * (datacol - upos[index]);

        index -= 264196;
    }
}


__attribute__((always_inline)) inline void forward_sweep_vec(index_t i,
    const index_t j,
    const index_t ishift,
    const index_t jshift,
    double *__restrict__ ccol,
    double *__restrict__ dcol,
    const double *__restrict__ wcon,
    const double *__restrict__ ustage,
    const double *__restrict__ upos,
    const double *__restrict__ utens,
    const double *__restrict__ utensstage) {

    vec_t ccol0, ccol1;
    vec_t dcol0, dcol1;
    vec_t ustage0, ustage1, ustage2;
    vec_t wcon0, wcon1;
    vec_t wcon_shift0, wcon_shift1;

    index_t index = i * 1 + j * 514;
    // k minimum
    {
        wcon_shift0 = loadu(&wcon[index + ishift * 1 + jshift * 514 + 264196]);
        wcon0 = load(&wcon[index + 264196]);
        vec_t gcv = double(0.25) * (wcon_shift0 + wcon0);
        vec_t cs = gcv * bet_m;

        ccol0 = gcv * bet_p;
        vec_t bcol = dtr_stage - ccol0;

        ustage0 = load(&ustage[index + 264196]);
        ustage1 = load(&ustage[index]);
        vec_t correction_term = -cs * (ustage0 - ustage1);
        dcol0 = dtr_stage * load(&upos[index]) + load(&utens[index]) + load(&utensstage[index]) + correction_term;

        vec_t divided = double(1.0) / bcol;
        ccol0 = ccol0 * divided;
        dcol0 = dcol0 * divided;

        store(&ccol[0], ccol0);
        store(&dcol[0], dcol0);

        index += 264196;
    }

    // k body
    for (index_t k = 1; k < 80 - 1; ++k) {
        

        ccol1 = ccol0;
        dcol1 = dcol0;
        ustage2 = ustage1;
        ustage1 = ustage0;
        wcon1 = wcon0;
        wcon_shift1 = wcon_shift0;

        vec_t gav = double(-0.25) * (wcon_shift1 + wcon1);
        wcon_shift0 = loadu(&wcon[index + ishift * 1 + jshift * 514 + 264196]);
        wcon0 = load(&wcon[index + 264196]);
        vec_t gcv = double(0.25) * (wcon_shift0 + wcon0);

        vec_t as = gav * bet_m;
        vec_t cs = gcv * bet_m;

        vec_t acol = gav * bet_p;
        ccol0 = gcv * bet_p;
        vec_t bcol = dtr_stage - acol - ccol0;

        ustage0 = load(&ustage[index + 264196]);
        vec_t correction_term = -as * (ustage2 - ustage1) - cs * (ustage0 - ustage1);
        dcol0 = dtr_stage * load(&upos[index]) + load(&utens[index]) + load(&utensstage[index]) + correction_term;

        vec_t divided = double(1.0) / (bcol - ccol1 * acol);
        ccol0 = ccol0 * divided;
        dcol0 = (dcol0 - dcol1 * acol) * divided;

        store(&ccol[k * 8], ccol0);
        store(&dcol[k * 8], dcol0);

        index += 264196;
    }

    // k maximum
    {
        ccol1 = ccol0;
        dcol1 = dcol0;
        ustage2 = ustage1;
        ustage1 = ustage0;
        wcon1 = wcon0;
        wcon_shift1 = wcon_shift0;

        vec_t gav = double(-0.25) * (wcon_shift1 + wcon1);

        vec_t as = gav * bet_m;

        vec_t acol = gav * bet_p;
        vec_t bcol = dtr_stage - acol;

        vec_t correction_term = -as * (ustage2 - ustage1);
        dcol0 = dtr_stage * load(&upos[index]) + load(&utens[index]) + load(&utensstage[index]) + correction_term;

        vec_t divided = double(1.0) / (bcol - ccol1 * acol);
        dcol0 = (dcol0 - dcol1 * acol) * divided;

        store(&ccol[79 * 8], ccol0);
        store(&dcol[79 * 8], dcol0);
    }
}


__attribute__((always_inline)) inline void backward_sweep_vec(index_t i,
    const index_t j,
    const double *__restrict__ ccol,
    const double *__restrict__ dcol,
    const double *__restrict__ upos,
    double *__restrict__ utensstage) {
    constexpr double dtr_stage = 3.0 / 20.0;

    vec_t datacol;

    index_t index = i * 1 + j * 514 + (80 - 1) * 264196;
    // k
    {
        datacol = load(&dcol[79 * 8]);
        store(&utensstage[index], dtr_stage * (datacol - load(&upos[index])));

        index -= 264196;
    }

    // k body
    for (index_t k = 80 - 2; k >= 0; --k) {
        datacol = load(&dcol[k * 8]) - load(&ccol[k * 8]) * datacol;
        store(&utensstage[index], dtr_stage * (datacol - load(&upos[index])));

        index -= 264196;
    }
}


void kernel_impl(
        double * __restrict__ ustage,
        double * __restrict__ upos,
        double * __restrict__ utens,
        double * __restrict__ utensstage,
        double * __restrict__ wcon,
        double * __restrict__ ccol,
        double * __restrict__ dcol,
        double * __restrict__ datacol
) {
    
#pragma omp parallel
    {
        alignas(0) double ccolb[640];
        alignas(0) double dcolb[640];

#pragma omp for collapse(2)
        for (index_t jb = 0; jb < 512; jb += 1) {
            for (index_t ib = 0; ib < 512; ib += 8) {
                    const index_t j = jb;
                    {
                        const index_t imax = std::min((index_t)512, ib + 8);

                        index_t i;
                        for (i = ib; i < imax - 7; i += 8) {
                            forward_sweep_vec(i, j, 1, 0, ccolb, dcolb, wcon, ustage, upos, utens, utensstage);
                            backward_sweep_vec(i, j, ccolb, dcolb, upos, utensstage);
                        }
                        for (; i < imax; ++i) {
                            forward_sweep(i, j, 1, 0, ccolb, dcolb, wcon, ustage, upos, utens, utensstage);
                            backward_sweep(i, j, ccolb, dcolb, upos, utensstage);
                        }
                    }
            }
        }
    }

}


extern "C" int kernel(
    double* time,
    long long* counter,
        double * __restrict__ ustage,
        double * __restrict__ upos,
        double * __restrict__ utens,
        double * __restrict__ utensstage,
        double * __restrict__ wcon,
        double * __restrict__ ccol,
        double * __restrict__ dcol,
        double * __restrict__ datacol
) {
    
    

    for (int dry_run = 0; dry_run < 0; ++dry_run) {
        kernel_impl(ustage, upos, utens, utensstage, wcon, ccol, dcol, datacol);
    }

    

    using clock = std::chrono::high_resolution_clock;
    auto start = clock::now();

    

    kernel_impl(ustage, upos, utens, utensstage, wcon, ccol, dcol, datacol);

    
    *counter = 0;
    

    auto stop = clock::now();
    *time = std::chrono::duration<double>(stop - start).count();
    return 0;
}
