/*
 * The chain latency probe (chain_probe.cuh) with the interval evaluation in
 * fixed point on the integer pipes (fixed_eval.cuh), beside elementwise.cu's
 * FP64 form: the two are bit-identical, and timing both on the same chains
 * shows which one a latency-bound kernel should use.
 */
#define MPRES_EVAL_FIXED_POINT 1
#include "kernels.h"
#include "mp_device.cuh"
#include "chain_probe.cuh"

MPRES_DEFINE_TABLES(probe_fx)

namespace mpres {
MPRES_CHAIN_PROBE_LAUNCHER(launch_chain_probe_fx)
} // namespace mpres
