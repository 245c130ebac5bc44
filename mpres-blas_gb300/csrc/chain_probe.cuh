/*
 * Latency probe of the reduction chains (mpres_probe_chain), included by
 * translation units that pick the interval evaluation with
 * MPRES_EVAL_FIXED_POINT: elementwise.cu (FP64, the form DOT, GEMV and SpMV
 * use) and probe_fx.cu (fixed point on the integer pipes, the form mp_gemm
 * uses), so both forms can be timed on the same chains.
 */
#ifndef MPRES_CHAIN_PROBE_CUH
#define MPRES_CHAIN_PROBE_CUH

namespace mpres {
namespace chainprobe {
using namespace dev;

/* the exponent mp_add gives x + y before any rounding (the expressions of
 * mp_add_common, src/arith/add.cuh:126-188); a rounding raises it by >= 1 */
template <int N> __device__ __forceinline__ int unrounded_sum_exp(const mp_t<N> &x, const mp_t<N> &y) {
    const Tables<N> &t = T<N>();
    int ex = x.exp, ey = y.exp;
    const int dexp = ex - ey;
    int gamma = dexp > 0 ? dexp : 0;
    int theta = dexp < 0 ? -dexp : 0;
    const int nzx = (!dnz(y.ev[1].frac) || (theta + y.ev[1].exp) < t.mp_j);
    const int nzy = (!dnz(x.ev[1].frac) || (gamma + x.ev[1].exp) < t.mp_j);
    gamma *= nzy;
    theta *= nzx;
    ex = (ex - gamma) * nzx;
    ey = (ey - theta) * nzy;
    return ex == 0 ? ey : ex;
}

/* Latency of the reduction chains, one warp alone on the GPU: lane l runs a
 * chain over elements l*len .. l*len+len-1 of
 *   kind 0: acc = acc + x*y   (mp_mul, mp_add: the DOT and GEMV step)
 *   kind 1: acc = acc + x     (mp_add alone: a step over precomputed products)
 *   kind 2: acc = acc + x*d   (mp_mul_d, mp_add: the SpMV step; y = double[])
 * Lane 0 writes the SM cycles of each step (clock64 between step ends; the next
 * step depends on the accumulator, so the deltas follow the dependent chain)
 * and how many lanes' product (bits 0-7) and sum (bits 8-15) rounded. */
template <int N>
__global__ void chain_probe(int kind, const void *x, const void *y, int len, long long *cycles, unsigned *rounds,
                            void *res) {
    const int lane = threadIdx.x;
    mp_t<N> acc;
    set_zero<N>(acc);
    long long prev = clock64();
    for (int t = 0; t < len; t++) {
        const long long i = (long long)lane * len + t;
        mp_t<N> a, p, s;
        load_aos<N>(a, x, i);
        bool pr = false;
        if (kind == 1) {
            p = a;
        } else if (kind == 0) {
            mp_t<N> b;
            load_aos<N>(b, y, i);
            mp_mul<N>(p, a, b);
            pr = p.exp != a.exp + b.exp;
        } else {
            const double d = __ldg(reinterpret_cast<const double *>(y) + i);
            const uint64_t u = dbits(d);
            const int dexp = dnz(d) ? (int)((u >> 52) & 2047) - 1075 : 0;
            mp_mul_d<N>(p, a, d);
            pr = p.exp != a.exp + dexp;
        }
        const int ue = unrounded_sum_exp<N>(acc, p);
        mp_add<N>(s, acc, p);
        const bool sr = s.exp != ue;
        acc = s;
        const unsigned np = __popc(__ballot_sync(0xffffffffu, pr)), ns = __popc(__ballot_sync(0xffffffffu, sr));
        const long long now = clock64();
        if (lane == 0) {
            cycles[t] = now - prev;
            rounds[t] = np | (ns << 8);
        }
        prev = clock64();
    }
    store_aos<N>(acc, res, lane);
}

/* Where a rounding's time goes, one warp alone: for `count` numbers per lane
 * (lane l takes digits of numbers l*count .. l*count+count-1, D[] the bits to
 * round away) lane 0 records per number the SM cycles of
 *   [0] rns_scale2pow(d, D), [1] rns_eval_compute_fast(d) (the rounding's two
 *   halves, mp_device.cuh's scale2pow and eval_fast), [2] one upward pairwise
 *   fraction sum psum_ru of the rounded residues, [3] the N modular products
 *   of one refinement step (s_i * RNS_POW2[k][i], k data dependent), and
 *   [4] rank_full of the input (the first scaling step's rank).
 * Results are written to `out` so nothing is optimised away. */
template <int N>
__global__ void round_parts_probe(const int *digits, const unsigned *D, int count, long long *cycles, int *out) {
    const Tables<N> &t = T<N>();
    const int lane = threadIdx.x;
    int acc = 0;
    for (int j = 0; j < count; j++) {
        const long long e = (long long)lane * count + j;
        int d[N], c[N];
#pragma unroll
        for (int i = 0; i < N; i++) d[i] = __ldg(digits + e * N + i);
        const unsigned bits = __ldg(D + e);
        __syncwarp();
        long long t0 = clock64();
#pragma unroll
        for (int i = 0; i < N; i++) c[i] = mulmod_i<N>(d[i], t.part_inv[i], i);
        const int rk = rank_full<N>(d, c);
        acc += rk;
        __syncwarp();
        long long t1 = clock64();
        scale2pow<N>(d, bits);
        acc += d[0];
        __syncwarp();
        long long t2 = clock64();
        er_t lo, up;
        eval_fast<N>(lo, up, d);
        acc += (int)up.exp;
        __syncwarp();
        long long t3 = clock64();
#pragma unroll
        for (int i = 0; i < N; i++) c[i] = mulmod_i<N>(d[i], t.part_inv[i], i);
        const double su = psum<N, true>([&](int i) { return __dmul_ru(u31_to_double((uint32_t)c[i]), t.recip_ru[i]); });
        acc += (int)(dbits(su) >> 40);
        __syncwarp();
        long long t4 = clock64();
        const int k = (int)(dbits(su) >> 52) & 63;
        const int *row = t.pow2 + (size_t)pow2_row_index<N>(k) * N;
#pragma unroll
        for (int i = 0; i < N; i++) c[i] = mulmod_i<N>(c[i], __ldg(row + i), i);
        acc += c[N - 1];
        __syncwarp();
        long long t5 = clock64();
        if (lane == 0) {
            cycles[j * 5 + 0] = t2 - t1;
            cycles[j * 5 + 1] = t3 - t2;
            cycles[j * 5 + 2] = t4 - t3;
            cycles[j * 5 + 3] = t5 - t4;
            cycles[j * 5 + 4] = t1 - t0;
        }
    }
    out[lane] = acc;
}

} // namespace chainprobe
} // namespace mpres

/* the host launchers of this translation unit's instantiations */
#define MPRES_ROUND_PROBE_LAUNCHER(NAME)                                                                      \
    cudaError_t NAME(int nmod, const int *digits, const unsigned *D, int count, long long *cycles, int *out,  \
                     cudaStream_t s) {                                                                        \
        switch (nmod) {                                                                                       \
        case 8: chainprobe::round_parts_probe<8><<<1, 32, 0, s>>>(digits, D, count, cycles, out); break;      \
        case 16: chainprobe::round_parts_probe<16><<<1, 32, 0, s>>>(digits, D, count, cycles, out); break;    \
        case 32: chainprobe::round_parts_probe<32><<<1, 32, 0, s>>>(digits, D, count, cycles, out); break;    \
        default: return cudaErrorInvalidValue;                                                                \
        }                                                                                                     \
        return cudaGetLastError();                                                                            \
    }
#define MPRES_CHAIN_PROBE_LAUNCHER(NAME)                                                                   \
    cudaError_t NAME(int nmod, int kind, const void *x, const void *y, int len, long long *cycles,         \
                     unsigned *rounds, void *res, cudaStream_t s) {                                        \
        switch (nmod) {                                                                                    \
        case 8: chainprobe::chain_probe<8><<<1, 32, 0, s>>>(kind, x, y, len, cycles, rounds, res); break;  \
        case 16: chainprobe::chain_probe<16><<<1, 32, 0, s>>>(kind, x, y, len, cycles, rounds, res); break; \
        case 32: chainprobe::chain_probe<32><<<1, 32, 0, s>>>(kind, x, y, len, cycles, rounds, res); break; \
        default: return cudaErrorInvalidValue;                                                             \
        }                                                                                                  \
        return cudaGetLastError();                                                                         \
    }

#endif
