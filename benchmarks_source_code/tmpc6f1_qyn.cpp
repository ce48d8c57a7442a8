

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
  using vec_t = double __attribute__((vector_size(1 * sizeof(double))));
  using ivec_t = index_t __attribute__((vector_size(1 * sizeof(index_t))));

  __attribute__((always_inline)) inline vec_t loadu(const double* ptr) {
#ifdef __clang__
    ptr = (double*)__builtin_assume_aligned(ptr, sizeof(double));
    vec_t v;
    for (int i = 0; i < 1; ++i)
      v[i] = ptr[i];
    return v;
#else
  using uvec_t = double __attribute__((vector_size(1 * sizeof(double)), aligned(sizeof(double))));
  return *(uvec_t*)ptr;
#endif
  }

  __attribute__((always_inline)) inline void storeu(double* ptr, vec_t v) {
#ifdef __clang__
    ptr = (double*)__builtin_assume_aligned(ptr, sizeof(double));
    for (int i = 0; i < 1; ++i)
      ptr[i] = v[i];
#else
    using uvec_t = double __attribute__((vector_size(1 * sizeof(double)), aligned(sizeof(double))));
    *(uvec_t*)ptr = v;
#endif
  }
    __attribute__((always_inline)) inline vec_t load(const double* ptr) { return loadu(ptr); }
    __attribute__((always_inline)) inline void store(double* ptr, vec_t v) { storeu(ptr, v); }
    __attribute__((always_inline)) inline void storent(double* ptr, vec_t v) { storeu(ptr, v); }

#ifdef __clang__
  __attribute__((always_inline)) inline vec_t select(ivec_t condition, vec_t v1, vec_t v2) {
    vec_t v;
    for (int i = 0; i < 1; ++i)
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
    
    constexpr index_t last = 1 * (512 - 1) +
                             516 * (512 - 1) +
                             266256 * (80 - 1);

    #pragma omp parallel for simd
    for (index_t index = 0; index <= last; ++index) {
        const auto inp_ij = inp[index];
                const auto inp_im1j = inp[index - 1];
                const auto inp_ip1j = inp[index + 1];
                const auto inp_ijm1 = inp[index - 516];
                const auto inp_ijp1 = inp[index + 516];
                const auto inp_im2j = inp[index - 2 * 1];
                const auto inp_im1jm1 = inp[index - 1 - 516];
                const auto inp_im1jp1 = inp[index - 1 + 516];
                const auto inp_ip2j = inp[index + 2 * 1];
                const auto inp_ip1jm1 = inp[index + 1 - 516];
                const auto inp_ip1jp1 = inp[index + 1 + 516];
                const auto inp_ijm2 = inp[index - 2 * 516];
                const auto inp_ijp2 = inp[index + 2 * 516];

                const auto lap_ij = 4 * inp_ij - inp_im1j
                                               - inp_ip1j
                                               - inp_ijm1
                                               - inp_ijp1;
                const auto lap_imj = 4 * inp_im1j - inp_im2j
                                                  - inp_ij
                                                  - inp_im1jm1
                                                  - inp_im1jp1;
                const auto lap_ipj = 4 * inp_ip1j - inp_ij
                                                  - inp_ip2j
                                                  - inp_ip1jm1
                                                  - inp_ip1jp1;
                const auto lap_ijm = 4 * inp_ijm1 - inp_im1jm1
                                                  - inp_ip1jm1
                                                  - inp_ijm2
                                                  - inp_ij;
                const auto lap_ijp = 4 * inp_ijp1 - inp_im1jp1
                                                  - inp_ip1jp1
                                                  - inp_ij
                                                  - inp_ijp2;

                auto flx_ij = lap_ipj - lap_ij;
                flx_ij = flx_ij * (inp_ip1j - inp_ij) > 0 ? 0 : flx_ij;

                auto flx_imj = lap_ij - lap_imj;
                flx_imj = flx_imj * (inp_ij - inp_im1j) > 0 ? 0 : flx_imj;

                auto fly_ij = lap_ijp - lap_ij;
                fly_ij = fly_ij * (inp_ijp1 - inp_ij) > 0 ? 0 : fly_ij;

                auto fly_ijm = lap_ij - lap_ijm;
                fly_ijm = fly_ijm * (inp_ij - inp_ijm1) > 0 ? 0 : fly_ijm;

                out[index] = inp_ij - coeff[index] * (flx_ij - flx_imj +
                                                      fly_ij - fly_ijm);
                
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
