/*
 * Conveyor entry points for the oracle build -- TEST INFRASTRUCTURE ONLY.
 * The conveyor library is not built for the oracle, so the three conveyor
 * variants report a set-up failure (-1.0), the reference's own convention
 * for "buffers could not be allocated" (apps/histo_src/histo_exstack.upc:58).
 */
#include <stdint.h>
#include "spmat.h"

double histo_conveyor(int64_t *pckindx, int64_t len, int64_t *lcounts) {
  (void)pckindx; (void)len; (void)lcounts; return -1.0;
}
double ig_conveyor(int64_t *tgt, int64_t *pckindx, int64_t l_num_req, int64_t *ltable) {
  (void)tgt; (void)pckindx; (void)l_num_req; (void)ltable; return -1.0;
}
double triangle_convey_push(int64_t *count, int64_t *sr, sparsemat_t *L, sparsemat_t *U, int64_t alg) {
  (void)count; (void)sr; (void)L; (void)U; (void)alg; return -1.0;
}
