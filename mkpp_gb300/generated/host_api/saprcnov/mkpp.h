/*
 * mkpp.h of the saprcnov library (libmkpp_saprcnov.so), generated from its plan.
 * The C ABI of include/mkpp.h plus the mechanism's sizes, as the header the
 * reference generates per mechanism defines them
 * (src/mkpp/templates/host_api/mkpp.h.j2:29-33).  A host model built against
 * that header puts this directory on its include path instead.
 */
#ifndef MKPP_GB300_SAPRCNOV_MKPP_H
#define MKPP_GB300_SAPRCNOV_MKPP_H

#include "../../../../include/mkpp.h"

#define MKPP_NUM_RATE_PARAMETERS 29
#define MKPP_NUM_SPECIES   96
#define MKPP_NUM_REACTIONS 187
#define MKPP_NUM_PHOTOLYSIS 29

/* Bytes of device memory that mkpp_gpu_integrate_noalloc's static scratch
 * holds on every GPU that loads this library, until the process exits. */
#define MKPP_NOALLOC_SCRATCH_BYTES (MKPP_NOALLOC_MAX_CELLS * 2111 * 8)

#endif
