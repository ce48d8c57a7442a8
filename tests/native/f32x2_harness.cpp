// Host build of the float-pair arithmetic (stencil_benchmarks_gb300/csrc/f32x2.cuh)
// for CPU tests: element-wise conversions and operations on double arrays.
#include "f32x2.cuh"

using sb::f32x2;

extern "C" {

void fx_split(const double* x, float* hi, float* lo, long n) {
    for (long q = 0; q < n; ++q) {
        const f32x2 v = sb::f32x2_from_double(x[q]);
        hi[q] = v.hi;
        lo[q] = v.lo;
    }
}

void fx_join(const float* hi, const float* lo, double* out, long n) {
    for (long q = 0; q < n; ++q) out[q] = sb::f32x2_to_double(f32x2(hi[q], lo[q]));
}

// op: 0 add, 1 sub, 2 mul, 3 div, 4 rcp(a), 5 cmp(a, b), 6 a * 4 (scale2<2>), 7 neg(a)
void fx_binop(int op, const double* a, const double* b, double* out, long n) {
    for (long q = 0; q < n; ++q) {
        const f32x2 x = sb::f32x2_from_double(a[q]), y = sb::f32x2_from_double(b[q]);
        f32x2 r(0);
        switch (op) {
            case 0: r = sb::add(x, y); break;
            case 1: r = sb::sub(x, y); break;
            case 2: r = sb::mul(x, y); break;
            case 3: r = sb::div(x, y); break;
            case 4: r = sb::rcp(x); break;
            case 5: out[q] = (double)sb::cmp(x, y); continue;
            case 6: r = sb::scale2<2>(x); break;
            case 7: r = -x; break;
        }
        out[q] = sb::f32x2_to_double(r);
    }
}

}  // extern "C"
