// Host build of the integer binary64 operations (stencil_benchmarks_gb300/
// csrc/softf64.cuh) for CPU tests: element-wise add / sub / mul / reciprocal
// on bit patterns, reporting whether the fast path took each case.
#include "softf64.cuh"

extern "C" {

// op: 0 add, 1 sub, 2 mul, 3 reciprocal of a (b unused).  taken[q] = 1 when
// the integer path produced out[q].
void sf_binop(int op, const uint64_t* a, const uint64_t* b, uint64_t* out, unsigned char* taken, long n) {
    for (long q = 0; q < n; ++q) {
        uint64_t r = 0;
        bool ok = false;
        switch (op) {
            case 0: ok = sb::sf::add(a[q], b[q], r); break;
            case 1: ok = sb::sf::sub(a[q], b[q], r); break;
            case 2: ok = sb::sf::mul(a[q], b[q], r); break;
            case 3: ok = sb::sf::rcp(a[q], r); break;
        }
        out[q] = r;
        taken[q] = ok ? 1 : 0;
    }
}

// ulps added to the reciprocal's float seed (the device's approximate
// reciprocal differs from the host's correctly rounded one by about 1 ulp)
void sf_set_rcp_perturb(int ulps) { sb::sf::rcp_seed_perturb() = ulps; }

}  // extern "C"
