/*
 * mkpp.h of the small_strato_rodas3 library (libmkpp_small_strato_rodas3.so), generated from its plan.
 * The C ABI of include/mkpp.h plus the mechanism's sizes, as the header the
 * reference generates per mechanism defines them
 * (src/mkpp/templates/host_api/mkpp.h.j2:29-33).  A host model built against
 * that header puts this directory on its include path instead.
 */
#ifndef MKPP_GB300_SMALL_STRATO_RODAS3_MKPP_H
#define MKPP_GB300_SMALL_STRATO_RODAS3_MKPP_H

#include "../../../../include/mkpp.h"

#define MKPP_NUM_RATE_PARAMETERS 4
#define MKPP_NUM_SPECIES   7
#define MKPP_NUM_REACTIONS 10
#define MKPP_NUM_PHOTOLYSIS 4

/* Bytes of device memory that mkpp_gpu_integrate_noalloc's static scratch
 * holds on every GPU that loads this library, until the process exits. */
#define MKPP_NOALLOC_SCRATCH_BYTES 8

#endif
