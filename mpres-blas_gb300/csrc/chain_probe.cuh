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

/* A leaf of the fraction sums, RU(s * recip_ru_i) (UP) or RD(s * recip_rd_i),
 * exactly, on the integer pipes: recip_i = R * 2^-83 with a 53-bit R, so the
 * product is the 84-bit integer P = s * R times 2^-83; rounding it to 53
 * significant bits (up: plus one unit when a dropped bit is set; down:
 * truncation) and assembling the double's fields gives the double that
 * __dmul_ru(s, recip_ru_i) / __dmul_rd(s, recip_rd_i) gives.  Measured as an
 * alternative to the FP64 leaves: the 64-bit integer products and the
 * normalisation cost more issue slots than the FP64 products they replace
 * (an 8-leaf upward sum took about 2480 cycles in context against 1250), so
 * the kernels keep __dmul_ru / __dmul_rd. */
template <int N, bool UP> __device__ __forceinline__ double int_leaf(uint32_t s, int i) {
    const Tables<N> &t = T<N>();
    const uint64_t R = UP ? t.recip_ru_m[i] : t.recip_rd_m[i];
    const uint64_t lo = (uint64_t)s * (uint32_t)R, hi = (uint64_t)s * (uint32_t)(R >> 32);
    const uint64_t plo = lo + (hi << 32);
    const uint64_t phi = (hi >> 32) + (plo < lo);
    if ((plo | phi) == 0) return 0.0;
    const int L = phi ? 128 - __clzll((long long)phi) : 64 - __clzll((long long)plo);
    uint64_t q;
    bool sticky;
    if (L > 53) {
        const int sh = L - 53; /* 1 .. 31 */
        q = (plo >> sh) | (phi << (64 - sh));
        sticky = (plo << (64 - sh)) != 0;
    } else {
        q = plo << (53 - L);
        sticky = false;
    }
    int e = L - 1 - 83; /* the value is in [2^e, 2^(e+1)) */
    if (UP && sticky) {
        q++;
        if (q >> 53) {
            q >>= 1;
            e++;
        }
    }
    return bdbl(((uint64_t)(e + 1023) << 52) | (q & ((1ull << 52) - 1)));
}

/* cycles of `reps` dependent fraction sums: form 0 = FP64 (the kernels' psum),
 * 1 = fixed point (fixed_eval.cuh), 2 = integer leaves and the FP64 tree */
template <int N>
__global__ void psum_probe(const int *digits, int form, int reps, long long *cycles, int *out) {
    const Tables<N> &t = T<N>();
    const int lane = threadIdx.x;
    int s[N];
#pragma unroll
    for (int i = 0; i < N; i++) s[i] = __ldg(digits + lane * N + i);
    int acc = 0;
    __syncwarp();
    const long long t0 = clock64();
    for (int r = 0; r < reps; r++) {
        uint64_t bits;
        if (form == 0) {
            bits = dbits(psum<N, true>([&](int i) { return __dmul_ru(u31_to_double((uint32_t)s[i]), t.recip_ru[i]); }));
        } else if (form == 1) {
            const fx f = fx_fraction_sum<N, true>(s);
            bits = f.lo ^ f.hi;
        } else {
            bits = dbits(psum<N, true>([&](int i) { return int_leaf<N, true>((uint32_t)s[i], i); }));
        }
#pragma unroll
        for (int i = 0; i < N; i++) s[i] ^= (int)((bits >> (i % 8)) & 1); /* every leaf of the next sum depends on this one */
        acc += (int)(bits >> 20);
    }
    const long long t1 = clock64();
    if (lane == 0) cycles[form] = (t1 - t0) / reps;
    out[lane] = acc + s[0];
}

/* int_leaf against __dmul_ru / __dmul_rd: out[4*i..] = {int RU, dmul RU, int RD, dmul RD} bits */
template <int N> __global__ void int_leaf_check(const int *digits, long long count, unsigned long long *out) {
    const Tables<N> &t = T<N>();
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count * N;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % N);
        const uint32_t s = (uint32_t)__ldg(digits + e);
        out[4 * e] = dbits(int_leaf<N, true>(s, i));
        out[4 * e + 1] = dbits(__dmul_ru(u31_to_double(s), t.recip_ru[i]));
        out[4 * e + 2] = dbits(int_leaf<N, false>(s, i));
        out[4 * e + 3] = dbits(__dmul_rd(u31_to_double(s), t.recip_rd[i]));
    }
}

/* the SM clock once v is computed: a shared-memory store of v (which waits for
 * it) and a block fence (which waits for the store) come first */
__device__ __forceinline__ long long clock_after(uint64_t v, volatile uint64_t *sink) {
    *sink = v;
    __threadfence_block();
    return clock64();
}

/* The phases of rns_eval_compute_fast (mp_device.cuh's eval_fast, FP64 form),
 * one warp alone, for `count` numbers per lane (lane l: digits of numbers
 * l*count .. l*count+count-1).  Lane 0 writes per number 4 + 3*12 counters:
 * [0] the part_inv products and the upward sum, [1] the number of refinement
 * steps, [2] the final downward sum, [3] the fence overhead of one clock_after;
 * then per refinement step j < 12: [4+3j] ceil(log2) and the row index, [5+3j]
 * the row load and the N modular products, [6+3j] the upward sum (leaves as
 * the library forms them, __dmul_ru). */
template <int N> __global__ void eval_phase_probe(const int *digits, int count, long long *cycles, int *out) {
    const Tables<N> &t = T<N>();
    __shared__ uint64_t sink[32];
    volatile uint64_t *mine = sink + threadIdx.x;
    const int lane = threadIdx.x;
    int acc = 0;
    for (int j = 0; j < count; j++) {
        long long c[4 + 36] = {};
        const long long e = (long long)lane * count + j;
        int s[N];
#pragma unroll
        for (int i = 0; i < N; i++) s[i] = __ldg(digits + e * N + i);
        long long t0 = clock_after((uint64_t)s[N - 1], mine);
        const long long t00 = clock_after((uint64_t)s[0], mine);
        c[3] = t00 - t0;
        t0 = t00;
#pragma unroll
        for (int i = 0; i < N; i++) s[i] = mulmod_i<N>(s[i], t.part_inv[i], i);
        double sumu = psum<N, true>([&](int i) { return __dmul_ru(u31_to_double((uint32_t)s[i]), t.recip_ru[i]); });
        sumu = d_frac<true>(sumu);
        long long t1 = clock_after(dbits(sumu), mine);
        c[0] = t1 - t0;
        int it = 0;
        for (int guard = 0; dbits(sumu) < dbits(t.eval_acc) && guard < 4096; guard++) {
            int k;
            if (!dnz(sumu)) {
                k = t.log2m;
            } else {
                const int cl = ceil_log2_d<N>(sumu);
                k = -(cl + 1) > t.ref_factor ? -(cl + 1) : t.ref_factor;
                k = pow2_row_index<N>(k < 0 ? 0 : k);
            }
            const long long ta = clock_after((uint64_t)k, mine);
            const int *row = t.pow2 + (size_t)k * N;
#pragma unroll
            for (int i = 0; i < N; i++) s[i] = mulmod_i<N>(s[i], __ldg(row + i), i);
            const long long tb = clock_after((uint64_t)s[N - 1] + (uint64_t)s[0], mine);
            sumu = psum<N, true>([&](int i) { return __dmul_ru(u31_to_double((uint32_t)s[i]), t.recip_ru[i]); });
            sumu = d_frac<true>(sumu);
            const long long tc = clock_after(dbits(sumu), mine);
            if (it < 12) {
                c[4 + 3 * it] = ta - t1;
                c[5 + 3 * it] = tb - ta;
                c[6 + 3 * it] = tc - tb;
            }
            t1 = tc;
            it++;
        }
        c[1] = it;
        const double suml =
            d_frac<false>(psum<N, false>([&](int i) { return __dmul_rd(u31_to_double((uint32_t)s[i]), t.recip_rd[i]); }));
        const long long t2 = clock_after(dbits(suml), mine);
        c[2] = t2 - t1;
        acc += (int)(dbits(suml) >> 33);
        if (lane == 0)
            for (int q = 0; q < 40; q++) cycles[(long long)j * 40 + q] = c[q];
    }
    out[lane] = acc;
}

} // namespace chainprobe
} // namespace mpres

/* the host launchers of this translation unit's instantiations */
#define MPRES_EVAL_PHASE_LAUNCHER(NAME)                                                                            \
    cudaError_t NAME(int nmod, const int *digits, int count, long long *cycles, int *out, cudaStream_t s) {     \
        switch (nmod) {                                                                                            \
        case 8: chainprobe::eval_phase_probe<8><<<1, 32, 0, s>>>(digits, count, cycles, out); break;               \
        case 16: chainprobe::eval_phase_probe<16><<<1, 32, 0, s>>>(digits, count, cycles, out); break;             \
        case 32: chainprobe::eval_phase_probe<32><<<1, 32, 0, s>>>(digits, count, cycles, out); break;             \
        default: return cudaErrorInvalidValue;                                                                     \
        }                                                                                                          \
        return cudaGetLastError();                                                                                 \
    }
#define MPRES_PSUM_PROBE_LAUNCHER(NAME)                                                                        \
    cudaError_t NAME(int nmod, int which, const int *digits, long long count, void *cycles_or_out, int *out,  \
                     cudaStream_t s) {                                                                          \
        if (which == 0) {                                                                                      \
            for (int f = 0; f < 3; f++) {                                                                      \
                if (nmod == 8) chainprobe::psum_probe<8><<<1, 32, 0, s>>>(digits, f, (int)count, (long long *)cycles_or_out, out); \
                else if (nmod == 16) chainprobe::psum_probe<16><<<1, 32, 0, s>>>(digits, f, (int)count, (long long *)cycles_or_out, out); \
                else if (nmod == 32) chainprobe::psum_probe<32><<<1, 32, 0, s>>>(digits, f, (int)count, (long long *)cycles_or_out, out); \
                else return cudaErrorInvalidValue;                                                             \
            }                                                                                                  \
            return cudaGetLastError();                                                                         \
        }                                                                                                      \
        const int g = 512;                                                                                     \
        if (nmod == 8) chainprobe::int_leaf_check<8><<<g, 256, 0, s>>>(digits, count, (unsigned long long *)cycles_or_out); \
        else if (nmod == 16) chainprobe::int_leaf_check<16><<<g, 256, 0, s>>>(digits, count, (unsigned long long *)cycles_or_out); \
        else if (nmod == 32) chainprobe::int_leaf_check<32><<<g, 256, 0, s>>>(digits, count, (unsigned long long *)cycles_or_out); \
        else return cudaErrorInvalidValue;                                                                     \
        return cudaGetLastError();                                                                             \
    }
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
