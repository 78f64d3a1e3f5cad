/* C-ABI wrapper around the reference's own host-compilable code
 * (TEST INFRASTRUCTURE ONLY; built by `make -C oracle ref` into oracle/_ref).
 * The reference's Thrust files (filter.cu, filter_by_mod.cu,
 * calc_mod_cands.cu, prepare_gen_mod.cu, gen_mod_pep.cu, prepare_scoring.cu,
 * sort.cu, prepare_ions_test.cu) are compiled unmodified from their own
 * sources with Thrust's CPP device system, so their extern "C" entry points
 * (algorithms.h:34-298) run on host memory.  This file only exposes the
 * inline combinatorics (combinatorics.h:59-134) and the C++-linkage
 * prepare_ions_test (prepare_ions_test.cu:47-55). */
#include <thrust/device_vector.h>
#include <cstdint>
#include <cstring>
#include "utils.h"
#include "algorithms.h"
#include "combinatorics.h"
#include "tests.h"

extern "C" uint32_t ref_choose(uint32_t n, uint32_t k) { return choose(n, k); }
extern "C" void ref_unrank_comb(uint32_t *ans, uint32_t n, uint32_t k, uint32_t rank) {
    unrankComb(ans, n, k, rank);
}
extern "C" void ref_prepare_ions(uint8_t *out, uint8_t *ions, uint32_t n, uint8_t *ma, uint32_t num_ma) {
    thrust::device_vector<uint8_t> r = prepare_ions_test(ions, n, ma, num_ma);
    thrust::copy(r.begin(), r.end(), out);
}
