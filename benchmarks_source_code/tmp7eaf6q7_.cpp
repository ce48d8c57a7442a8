

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




void kernel_impl(
        double * __restrict__ inp,
        double * __restrict__ coeff,
        double * __restrict__ out
) {
    
#pragma omp parallel for collapse(3)
  for (index_t kb = 0; kb < 80; kb += 1) {
    for (index_t jb = 0; jb < 512; jb += 8) {
      for (index_t ib = 0; ib < 512; ib += 8) {
          const index_t imax = std::min(512 - ib, (index_t)8);
          const index_t jmax = std::min(512 - jb, (index_t)8);
          const index_t k = 0;
          {

            for (index_t j = 0; j < jmax; ++j) {
              constexpr vec_t zero_vec = { 0, 0, 0, 0, 0, 0, 0, 0 };
              index_t i;
              for (i = 0; i < imax - 7; i += 8) {
                const index_t index = (ib + i) * 1 + (jb + j) * 516 + (kb + k) * 266256;

                const vec_t inp_ij = load(&inp[index]);
                const vec_t inp_im1j = loadu(&inp[index - 1]);
                const vec_t inp_ip1j = loadu(&inp[index + 1]);
                const vec_t inp_ijm1 = load(&inp[index - 516]);
                const vec_t inp_ijp1 = load(&inp[index + 516]);
                const vec_t inp_im2j = loadu(&inp[index - 2 * 1]);
                const vec_t inp_im1jm1 = loadu(&inp[index - 1 - 516]);
                const vec_t inp_im1jp1 = loadu(&inp[index - 1 + 516]);
                const vec_t inp_ip2j = loadu(&inp[index + 2 * 1]);
                const vec_t inp_ip1jm1 = loadu(&inp[index + 1 - 516]);
                const vec_t inp_ip1jp1 = loadu(&inp[index + 1 + 516]);
                const vec_t inp_ijm2 = load(&inp[index - 2 * 516]);
                const vec_t inp_ijp2 = load(&inp[index + 2 * 516]);

                const vec_t lap_ij = 4 * inp_ij - inp_im1j - inp_ip1j -
                inp_ijm1 - inp_ijp1;
                const vec_t lap_imj = 4 * inp_im1j - inp_im2j -
                    inp_ij - inp_im1jm1 -
                    inp_im1jp1;
                const vec_t lap_ipj = 4 * inp_ip1j - inp_ij -
                    inp_ip2j - inp_ip1jm1 -
                    inp_ip1jp1;
                const vec_t lap_ijm = 4 * inp_ijm1 - inp_im1jm1 -
                    inp_ip1jm1 - inp_ijm2 -
                    inp_ij;
                const vec_t lap_ijp = 4 * inp_ijp1 - inp_im1jp1 -
                    inp_ip1jp1 - inp_ij -
                    inp_ijp2;

                vec_t flx_ij = lap_ipj - lap_ij;
                flx_ij = select(flx_ij * (inp_ip1j - inp_ij) > 0, zero_vec, flx_ij);

                vec_t flx_imj = lap_ij - lap_imj;
                flx_imj = select(flx_imj * (inp_ij - inp_im1j) > 0, zero_vec, flx_imj);

                vec_t fly_ij = lap_ijp - lap_ij;
                fly_ij = select(fly_ij * (inp_ijp1 - inp_ij) > 0, zero_vec, fly_ij);

                vec_t fly_ijm = lap_ij - lap_ijm;
                fly_ijm = select(fly_ijm * (inp_ij - inp_ijm1) > 0, zero_vec, fly_ijm);

                vec_t out_ij = inp_ij - load(&coeff[index]) * (flx_ij - flx_imj +
                                                               fly_ij - fly_ijm);
                storent(&out[index], out_ij);
              }

              for (; i < imax; ++i) {
                const index_t index = (ib + i) * 1 + (jb + j) * 516 + (kb + k) * 266256;

                const double inp_ij = inp[index];
                const double inp_im1j = inp[index - 1];
                const double inp_ip1j = inp[index + 1];
                const double inp_ijm1 = inp[index - 516];
                const double inp_ijp1 = inp[index + 516];
                const double inp_im2j = inp[index - 2 * 1];
                const double inp_im1jm1 = inp[index - 1 - 516];
                const double inp_im1jp1 = inp[index - 1 + 516];
                const double inp_ip2j = inp[index + 2 * 1];
                const double inp_ip1jm1 = inp[index + 1 - 516];
                const double inp_ip1jp1 = inp[index + 1 + 516];
                const double inp_ijm2 = inp[index - 2 * 516];
                const double inp_ijp2 = inp[index + 2 * 516];

                const double lap_ij = 4 * inp_ij - inp_im1j - inp_ip1j -
                inp_ijm1 - inp_ijp1;
                const double lap_imj = 4 * inp_im1j - inp_im2j -
                    inp_ij - inp_im1jm1 -
                    inp_im1jp1;
                const double lap_ipj = 4 * inp_ip1j - inp_ij -
                    inp_ip2j - inp_ip1jm1 -
                    inp_ip1jp1;
                const double lap_ijm = 4 * inp_ijm1 - inp_im1jm1 -
                    inp_ip1jm1 - inp_ijm2 -
                    inp_ij;
                const double lap_ijp = 4 * inp_ijp1 - inp_im1jp1 -
                    inp_ip1jp1 - inp_ij -
                    inp_ijp2;

                double flx_ij = lap_ipj - lap_ij;
                flx_ij = flx_ij * (inp_ip1j - inp_ij) > 0 ? 0 : flx_ij;

                double flx_imj = lap_ij - lap_imj;
                flx_imj = flx_imj * (inp_ij - inp_im1j) > 0 ? 0 : flx_imj;

                double fly_ij = lap_ijp - lap_ij;
                fly_ij = fly_ij * (inp_ijp1 - inp_ij) > 0 ? 0 : fly_ij;

                double fly_ijm = lap_ij - lap_ijm;
                fly_ijm = fly_ijm * (inp_ij - inp_ijm1) > 0 ? 0 : fly_ijm;

                out[index] = inp_ij - coeff[index] * (flx_ij - flx_imj +
                                        fly_ij - fly_ijm);
              }
              /* nonsense data modification to avoid break in access stream and thus hardware prefetching failure */
              if (ib + 8 >= 512) {
                const index_t index = (ib + imax) * 1 + (jb + j) * 516 + (kb + k) * 266256;
                out[index] = inp[index] + inp[index + 1032] + coeff[index];
              }
            }
          }
      }
    }
  }

}


extern "C" int kernel(
    double* time,
    long long* counter,
        double * __restrict__ inp,
        double * __restrict__ coeff,
        double * __restrict__ out
) {
    
    

    for (int dry_run = 0; dry_run < 0; ++dry_run) {
        kernel_impl(inp, coeff, out);
    }

    

    using clock = std::chrono::high_resolution_clock;
    auto start = clock::now();

    

    kernel_impl(inp, coeff, out);

    
    *counter = 0;
    

    auto stop = clock::now();
    *time = std::chrono::duration<double>(stop - start).count();
    return 0;
}
