/*
 * Diagnostic entry points of libmpres_gb300.so (no counterpart in the
 * reference, which has no benchmarking API).  They launch throughput
 * microkernels on `stream` and return at once; the caller times them with
 * events.  Each thread performs 8 independent chains of `iters` operations:
 *   mpres_probe_mulmod: blocks*threads*iters*8 Barrett modular products
 *                       (the residue reduction every RNS kernel uses);
 *   mpres_probe_dadd:   blocks*threads*iters*8 directed-rounding double adds.
 * `sink` is a device buffer of at least 8 bytes that the kernels may write.
 */
#ifndef MPRES_GB300_PROBE_H
#define MPRES_GB300_PROBE_H

#include <stddef.h>

#include "mpres_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

int mpres_probe_mulmod(int blocks, int threads, long long iters, void *sink, void *stream);
int mpres_probe_dadd(int blocks, int threads, long long iters, void *sink, void *stream);
/* Latency of one dependent operation in SM cycles, measured by one thread over
 * `iters` operations: which 0 = __dadd_rd, 1 = Barrett modular product,
 * 2 = 64-bit shift-add; out = device double[2], out[0] receives the cycles. */
int mpres_probe_latency(int which, long long iters, void *out, void *stream);

/* out[i] = ceil(log2(x[i])) with the CUDA math library, the expression the
 * reference's interval-evaluation refinement loop evaluates on the device
 * (src/rns.cuh:848, :913); x and out are double[count] in device memory. */
int mpres_probe_ceil_log2(const double *x, double *out, size_t count, void *stream);

/* Self-checks of the exact replacements the kernels use for CUDA operations
 * (each writes the replacement's result next to the CUDA operation's):
 *   which 0: directed division by the set's RNS_EVAL_UNIT bounds, a = double[count],
 *            out = double[4*count]: {div_rd, __ddiv_rd, div_ru, __ddiv_ru};
 *   which 1: exponent-field scaling, a = double[count], b = int[count],
 *            out = double[2*count]: {scale2(a, b), scalbn(a, b)};
 *   which 2: ceil(log2) of fixed-point fractions, a = double[count] (multiples of
 *            2^-83 below 1), out = int[2*count]: {from bits, ceil(log2(a))};
 *   which 3: ceil(log2) of any positive doubles, a = double[count],
 *            out = int[2*count]: {from bits, ceil(log2(a))}.
 * All pointers are device memory. */
int mpres_probe_check(int which, int nmod, const void *a, const void *b, void *out, size_t count, void *stream);

/* Latency of the reduction chains on one warp running alone: 32 chains of len
 * steps, lane l over elements l*len .. l*len+len-1 of
 *   kind 0: acc = acc + x[i]*y[i]   (cuda::mp_mul + cuda::mp_add, the DOT/GEMV step)
 *   kind 1: acc = acc + x[i]        (cuda::mp_add alone)
 *   kind 2: acc = acc + x[i]*y[i]   (cuda::mp_mul_d + cuda::mp_add, the SpMV step; y = double[])
 * x, y: AoS mp_float_t[32*len] (y double[32*len] for kind 2); cycles: long long[len]
 * receives the SM cycles of each step; rounds: unsigned[len] the number of lanes
 * whose product (bits 0-7) and sum (bits 8-15) rounded at that step; result:
 * mp_float_t[32], each lane's sum.  All pointers are device memory.
 * kind + MPRES_PROBE_FIXED_POINT runs the same chains with the interval
 * evaluation in fixed point on the integer pipes instead of FP64 (same bits). */
#define MPRES_PROBE_FIXED_POINT 16
int mpres_probe_chain(int nmod, int kind, const void *x, const void *y, int len, long long *cycles,
                      unsigned *rounds, void *result, void *stream);

/* Where the time of a rounding goes, one warp alone: digits = int[32*count*nmod]
 * (lane l takes numbers l*count .. l*count+count-1), D = unsigned[32*count]
 * bits to round away; cycles = long long[count*5] receives lane 0's SM cycles
 * per number of {rns_scale2pow, rns_eval_compute_fast, one upward fraction
 * sum, the modular products of one refinement step, rank_full}; out = int[32]
 * (a checksum).  Device memory. */
int mpres_probe_rounding(int nmod, const int *digits, const unsigned *D, int count, long long *cycles, int *out,
                         void *stream);

/* The upward fraction sum of the interval evaluation three ways, exact and
 * bit-identical: which 0 times `count` dependent sums on one warp for each form
 * (digits = int[32*nmod] residues, result = long long[3] cycles per sum of
 * {FP64 as the reference, fixed point, integer leaves + FP64 tree}, out =
 * int[32] checksum); which 1 checks the integer leaves against __dmul_ru /
 * __dmul_rd on digits = int[count*nmod], result = unsigned long long[4*count*nmod]
 * {integer RU, __dmul_ru, integer RD, __dmul_rd} bits.  Device memory. */
int mpres_probe_fraction_sum(int nmod, int which, const int *digits, long long count, void *result, int *out,
                             void *stream);

/* The phases of the interval evaluation rns_eval_compute_fast, one warp alone:
 * digits = int[32*count*nmod] (lane l takes numbers l*count ..
 * l*count+count-1); cycles = long long[40*count] receives lane 0's SM cycles
 * per number: {initial products and upward sum, refinement steps taken, final
 * downward sum, clock-fence overhead, then for each of up to 12 refinement
 * steps: ceil(log2) and row index, row load and modular products, upward
 * sum}; out = int[32] checksum.  Device memory. */
int mpres_probe_eval_phases(int nmod, const int *digits, int count, long long *cycles, int *out, void *stream);

/* mp_gemm (no transposes, 32 moduli) in its split form with an event between
 * its phases: ms = float[7] receives the time of each -- W(A), W(B), their limb
 * planes, the scalar chain, the modular product on the tensor cores, the
 * epilogue, the per-output chain of the outputs that leave that form -- after
 * the call has completed on `stream`.  Same arguments and results as mpres_gemm
 * otherwise. */
int mpres_probe_gemm_phases(int nmod, int m, int n, int k, const mp_array_t *alpha, const mp_array_t *A, int lda,
                            const mp_array_t *B, int ldb, const mp_array_t *beta, mp_array_t *C, int ldc, float *ms,
                            void *stream);

/* Element-wise device arithmetic over AoS mp_float_t vectors (device memory), one
 * element per thread: the device functions the BLAS kernels are built from,
 * exposed so that each can be checked against the reference on its own.
 *   MPRES_OP_ADD:   r[i] = x[i] + y[i]   cuda::mp_add (src/arith/add.cuh:190-202)
 *   MPRES_OP_MUL:   r[i] = x[i] * y[i]   cuda::mp_mul (src/arith/mul.cuh:71-80)
 *   MPRES_OP_MUL_D: r[i] = x[i] * d[i]   cuda::mp_mul_d (src/arith/muld.cuh:59-74), y = double[count] */
#define MPRES_OP_ADD 0
#define MPRES_OP_MUL 1
#define MPRES_OP_MUL_D 2
int mpres_elementwise(int nmod, int op, const void *x, const void *y, void *r, size_t count, void *stream);

/* cuda::rns_scale2pow (src/rns.cuh:1132-1158): out = digits / 2^D[i], digits and out
 * int[count * nmod] in device memory. */
int mpres_rns_scale2pow(int nmod, const int *digits, const unsigned *D, int *out, size_t count, void *stream);

/* cuda::rns_eval_compute (fast = 0, src/rns.cuh:797-868) or rns_eval_compute_fast
 * (fast = 1, :878-933): interval evaluation of digits[count * nmod] into low[count],
 * upp[count] (er_float_t, device memory). */
int mpres_rns_eval(int nmod, int fast, const int *digits, void *low, void *upp, size_t count, void *stream);

#ifdef __cplusplus
}
#endif

#endif
