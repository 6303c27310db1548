// ===========================================================================
// Standalone build of the synthetic-data generator -- MEASUREMENT
// INFRASTRUCTURE ONLY.
//
// bench.py's CPU arms (the reference arm and the cpu_baseline leg) draw their
// input from the BUSseq generative model like the GPU arm does, but must not
// map the product library (libbusseq_gb300.so) while they run: their process
// is meant to hold only the checker side.  This file compiles the product's
// generator source (busseq_gpu_gb300/csrc/simulate.cpp, host code only) into
// oracle/lib/libsim.so together with the one library function it calls, so the
// same seed gives the same counts in both libraries
// (tests/test_bench_baselines.py checks that).
// ===========================================================================
#include <stdio.h>
#include <string.h>

static char g_err[512];

extern "C" int busseq_internal_set_error(int code, const char* msg) {
  snprintf(g_err, sizeof g_err, "%s", msg ? msg : "");
  return code;
}

extern "C" const char* sim_last_error() { return g_err; }

#include "simulate.cpp"
