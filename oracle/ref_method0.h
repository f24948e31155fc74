/* Forced-include header for compiling the reference's tc/bs_tc/bs_tc.cu, unmodified, with
 * its method 0 (ListIntersectionKernel, bs_tc.cu:120-148) instead of the method 1 its
 * shipped tc/rt_tc/include/config.h selects. config.h is included here first; its
 * `#pragma once` makes the source's own include of it a no-op, and the method is redefined.
 * TEST INFRASTRUCTURE ONLY (the reference's GPU kernel as a same-box data point). */
#include "config.h"
#undef RTTC_METHOD
#define RTTC_METHOD 0
