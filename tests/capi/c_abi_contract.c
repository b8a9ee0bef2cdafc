/* The reference's C-ABI contract tests (tests/contract/test_c_abi.cpp:9-80:
 * handle lifecycle and error handling, state binding validation, batch
 * photolysis binding) as a C11 program built against a mechanism's generated
 * mkpp.h and linked to its library (TEST INFRASTRUCTURE ONLY; run by
 * tests/test_capi_contract.py).  No call here computes, so no GPU is needed.
 * Prints "ok" and exits 0 when every expectation holds. */
#include <stdio.h>
#include <stdlib.h>

#include "mkpp.h"

#define EXPECT(c)                                                 \
  do {                                                            \
    if (!(c)) {                                                   \
      fprintf(stderr, "%s:%d: expected %s\n", __FILE__, __LINE__, #c); \
      return 1;                                                   \
    }                                                             \
  } while (0)

static double* filled(size_t n, double v) {
  double* p = (double*)malloc(n * sizeof(double));
  for (size_t i = 0; i < n; ++i) p[i] = v;
  return p;
}

static int lifecycle(void) {
  mkpp_handle_t h = NULL;
  EXPECT(mkpp_initialize(h) == MKPP_ERROR_NULL_POINTER);
  EXPECT(mkpp_create_handle(&h, 10) == MKPP_SUCCESS);
  EXPECT(h != NULL);
  EXPECT(mkpp_initialize(h) == MKPP_SUCCESS);
  size_t count = 0;
  EXPECT(mkpp_get_species_count(h, &count) == MKPP_SUCCESS && count == (size_t)MKPP_NUM_SPECIES);
  EXPECT(mkpp_get_reaction_count(h, &count) == MKPP_SUCCESS && count == (size_t)MKPP_NUM_REACTIONS);
  EXPECT(mkpp_get_photolysis_count(h, &count) == MKPP_SUCCESS && count == (size_t)MKPP_NUM_PHOTOLYSIS);
  EXPECT(mkpp_destroy_handle(h) == MKPP_SUCCESS);
  return 0;
}

static int state_binding(void) {
  const size_t cells = 5, ns = MKPP_NUM_SPECIES;
  mkpp_handle_t h = NULL;
  EXPECT(mkpp_create_handle(&h, cells) == MKPP_SUCCESS);
  EXPECT(mkpp_initialize(h) == MKPP_SUCCESS);
  double *conc = filled(cells * ns, 1.0e-9), *temp = filled(cells, 298.15), *pres = filled(cells, 101325.0),
         *rho = filled(cells, 2.45e19);
  EXPECT(mkpp_set_state_ptrs(h, NULL, temp, pres, rho) == MKPP_ERROR_NULL_POINTER);
  EXPECT(mkpp_set_state_ptrs(h, conc, temp, pres, rho) == MKPP_SUCCESS);
  EXPECT(mkpp_destroy_handle(h) == MKPP_SUCCESS);
  free(conc), free(temp), free(pres), free(rho);
  return 0;
}

static int photolysis_binding(void) {
  const size_t cells = 100, ns = MKPP_NUM_SPECIES;
  const size_t nph = MKPP_NUM_PHOTOLYSIS > 0 ? MKPP_NUM_PHOTOLYSIS : 1;
  mkpp_handle_t h = NULL;
  EXPECT(mkpp_create_handle(&h, cells) == MKPP_SUCCESS);
  EXPECT(mkpp_initialize(h) == MKPP_SUCCESS);
  double *conc = filled(cells * ns, 1.0e-9), *temp = filled(cells, 298.15), *pres = filled(cells, 101325.0),
         *rho = filled(cells, 2.45e19), *photo = filled(cells * nph, 1.0e-5), *rh = filled(cells, 70.0),
         *sa = filled(cells, 1.0e-4);
  EXPECT(mkpp_set_state_ptrs(h, conc, temp, pres, rho) == MKPP_SUCCESS);
  /* As in the reference (mkpp_c_api.cpp.j2:207-210): photolysis rates alone
   * bind only when they are the whole runtime parameter array. */
  if (MKPP_NUM_RATE_PARAMETERS > MKPP_NUM_PHOTOLYSIS) {
    EXPECT(mkpp_set_photolysis_ptrs(h, photo) == MKPP_ERROR_INVALID_ARGUMENT);
  } else {
    EXPECT(mkpp_set_photolysis_ptrs(h, photo) == MKPP_SUCCESS);
  }
  EXPECT(mkpp_set_aerosol_ptrs(h, rh, sa) == MKPP_SUCCESS);
  EXPECT(mkpp_destroy_handle(h) == MKPP_SUCCESS);
  free(conc), free(temp), free(pres), free(rho), free(photo), free(rh), free(sa);
  return 0;
}

int main(void) {
  if (lifecycle() || state_binding() || photolysis_binding()) return 1;
  puts("ok");
  return 0;
}
