// Host build of the integer binary64 operations (stencil_benchmarks_gb300/
// csrc/softf64.cuh) for CPU tests: element-wise add / sub / mul on bit
// patterns, reporting whether the fast path took each case.
#include "softf64.cuh"

extern "C" {

// op: 0 add, 1 sub, 2 mul.  taken[q] = 1 when the integer path produced out[q].
void sf_binop(int op, const uint64_t* a, const uint64_t* b, uint64_t* out, unsigned char* taken, long n) {
    for (long q = 0; q < n; ++q) {
        uint64_t r = 0;
        bool ok = false;
        switch (op) {
            case 0: ok = sb::sf::add(a[q], b[q], r); break;
            case 1: ok = sb::sf::sub(a[q], b[q], r); break;
            case 2: ok = sb::sf::mul(a[q], b[q], r); break;
        }
        out[q] = r;
        taken[q] = ok ? 1 : 0;
    }
}

}  // extern "C"
