// flop_count.cpp -- TEST INFRASTRUCTURE ONLY: the counters of the op-counting
// build of the oracle (see flop_count.h) and their C entry point.
#include "flop_count.h"

unsigned long long g_oracle_ops[OC_N];

// Copy the counters (add/subtract, multiply, divide, sqrt, compare, min/max,
// abs) into out[7]; with reset, zero them afterwards.
extern "C" void oracle_op_counts(unsigned long long* out, int reset) {
  for (int k = 0; k < OC_N; k++) {
    if (out) out[k] = g_oracle_ops[k];
    if (reset) g_oracle_ops[k] = 0;
  }
}
