/*
 * Host-side stand-ins for the CUDA language features used by the reference
 * library's device code, so that its unmodified headers compile with g++ and
 * its device functions and kernels run on the CPU:
 *
 *   - execution-space qualifiers become no-ops (`__shared__` arrays declared
 *     `extern` resolve to one block-wide global array defined by the harness);
 *   - threadIdx/blockIdx/blockDim/gridDim are globals set by a launcher that
 *     runs every thread of a block as a ucontext coroutine, so __syncthreads()
 *     is a real block-wide barrier;
 *   - the directed-rounding intrinsics (__dadd_rd, __dmul_ru, __ddiv_rd, ...)
 *     are IEEE-754 operations performed under fesetround(), which is exactly
 *     what the CUDA intrinsics specify;
 *   - the memory API (cudaMalloc, cudaMemcpy, cudaMemcpyToSymbol) is host
 *     memory.
 *
 * Test infrastructure only: it builds the reference under oracle/_ref/ to pin
 * the oracle; nothing in the product links it.
 */
#ifndef ORACLE_CUDA_EMU_H
#define ORACLE_CUDA_EMU_H

#include <cfenv>
#include <cstdint>
#include <iostream>
#include <string>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <ucontext.h>
#include <vector>

#define __host__
#define __device__
#define __global__
#define __constant__
#define __shared__
#define __forceinline__ inline
#define __noinline__

struct int4 { int x, y, z, w; };
struct uint3 { unsigned int x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};

extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
                      cudaMemcpyDeviceToDevice };
enum cudaFuncCache { cudaFuncCachePreferNone, cudaFuncCachePreferShared };
inline const char *cudaGetErrorString(cudaError_t) { return "no error"; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaDeviceReset() { return cudaSuccess; }
template <class T> inline cudaError_t cudaMalloc(T **p, size_t sz) { *p = (T *)calloc(1, sz ? sz : 1); return 0; }
inline cudaError_t cudaFree(void *p) { free(p); return 0; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t sz, cudaMemcpyKind) { memcpy(d, s, sz); return 0; }
template <class S, class T> inline cudaError_t cudaMemcpyToSymbol(S &sym, const T *src, size_t sz) {
    memcpy((void *)&sym, (const void *)src, sz);
    return 0;
}
template <class F> inline cudaError_t cudaFuncSetCacheConfig(F, cudaFuncCache) { return 0; }

/* ---- directed rounding: IEEE operations under an explicit rounding mode ---- */
#define ORACLE_DIRECTED(name, op, mode)                                   \
    static inline double name(double a, double b) {                       \
        volatile double va = a, vb = b;                                   \
        fesetround(mode);                                                 \
        volatile double r = va op vb;                                     \
        fesetround(FE_TONEAREST);                                         \
        return r;                                                         \
    }
ORACLE_DIRECTED(__dadd_rd, +, FE_DOWNWARD)
ORACLE_DIRECTED(__dadd_ru, +, FE_UPWARD)
ORACLE_DIRECTED(__dadd_rn, +, FE_TONEAREST)
ORACLE_DIRECTED(__dsub_rd, -, FE_DOWNWARD)
ORACLE_DIRECTED(__dsub_ru, -, FE_UPWARD)
ORACLE_DIRECTED(__dmul_rd, *, FE_DOWNWARD)
ORACLE_DIRECTED(__dmul_ru, *, FE_UPWARD)
ORACLE_DIRECTED(__dmul_rn, *, FE_TONEAREST)
ORACLE_DIRECTED(__ddiv_rd, /, FE_DOWNWARD)
ORACLE_DIRECTED(__ddiv_ru, /, FE_UPWARD)
#undef ORACLE_DIRECTED

/* ---- CUDA's log2 as the device code sees it ----
 * The reference's device code uses log2 only for ceil(log2(sumu)) in its
 * interval-evaluation refinement loop (src/rns.cuh:848, :913).  CUDA's log2 can
 * be one ulp off the exact value within a few ulps of a power of two, which
 * changes that ceiling; cuda_log2_table.h lists those deviations as measured on
 * the GPU.  Unqualified calls inside namespace cuda resolve to this function,
 * which returns a value whose ceiling is CUDA's; host code keeps the C library's. */
#include "cuda_log2_table.h"
namespace emu_log2 {
    inline int delta(int e, long long steps) {
        for (int r = 0; r < ORA_CUDA_LOG2_RUNS; r++)
            if (ORA_CUDA_LOG2_TABLE[r][0] == e && steps >= ORA_CUDA_LOG2_TABLE[r][1] &&
                steps <= ORA_CUDA_LOG2_TABLE[r][2])
                return ORA_CUDA_LOG2_TABLE[r][3];
        return 0;
    }
    inline long long bits(double d) { long long u; memcpy(&u, &d, 8); return u; }
}
namespace cuda {
    inline double log2(double x) {
        int e;
        double m = frexp(x, &e);
        double exact = (m == 0.5) ? e - 1 : e;
        e -= 1;
        int d = emu_log2::delta(e, emu_log2::bits(x) - emu_log2::bits(ldexp(1.0, e)));
        if (!d) d = emu_log2::delta(e + 1, emu_log2::bits(x) - emu_log2::bits(ldexp(1.0, e + 1)));
        return exact + d - 0.5;
    }
}

/* ---- block execution: one coroutine per thread, __syncthreads() yields ---- */
namespace emu {
    struct Block {
        std::vector<ucontext_t> ctx;
        std::vector<char> done;
        std::vector<uint3> tid;
        ucontext_t sched;
        int cur = -1;
        std::function<void()> body;
    };
    extern Block *g_block;
    extern std::vector<char> g_stacks;
    constexpr size_t kStack = 256 * 1024;

    inline void trampoline() {
        Block *b = g_block;
        b->body();
        b->done[b->cur] = 1;
        swapcontext(&b->ctx[b->cur], &b->sched);
    }

    /* Runs body for every thread of every block of the grid. */
    inline void launch(dim3 grid, dim3 block, const std::function<void()> &body, bool barriers) {
        gridDim = grid;
        blockDim = block;
        const int nt = block.x * block.y * block.z;
        for (unsigned bz = 0; bz < grid.z; bz++)
        for (unsigned by = 0; by < grid.y; by++)
        for (unsigned bx = 0; bx < grid.x; bx++) {
            blockIdx = {bx, by, bz};
            if (!barriers) {
                for (int t = 0; t < nt; t++) {
                    threadIdx = {(unsigned)(t % block.x), (unsigned)((t / block.x) % block.y),
                                 (unsigned)(t / (block.x * block.y))};
                    body();
                }
                continue;
            }
            Block b;
            b.ctx.resize(nt);
            b.done.assign(nt, 0);
            b.tid.resize(nt);
            b.body = body;
            if (g_stacks.size() < nt * kStack) g_stacks.resize(nt * kStack);
            g_block = &b;
            for (int t = 0; t < nt; t++) {
                b.tid[t] = {(unsigned)(t % block.x), (unsigned)((t / block.x) % block.y),
                            (unsigned)(t / (block.x * block.y))};
                getcontext(&b.ctx[t]);
                b.ctx[t].uc_stack.ss_sp = &g_stacks[t * kStack];
                b.ctx[t].uc_stack.ss_size = kStack;
                b.ctx[t].uc_link = nullptr;
                makecontext(&b.ctx[t], (void (*)())trampoline, 0);
            }
            bool all_done = false;
            while (!all_done) {
                all_done = true;
                for (int t = 0; t < nt; t++) {
                    if (b.done[t]) continue;
                    b.cur = t;
                    threadIdx = b.tid[t];
                    swapcontext(&b.sched, &b.ctx[t]);
                    if (!b.done[t]) all_done = false;
                }
            }
            g_block = nullptr;
        }
    }
}

inline void __syncthreads() {
    emu::Block *b = emu::g_block;
    if (!b) return; /* barrier-free launch: nothing to wait for */
    swapcontext(&b->ctx[b->cur], &b->sched);
}

#endif
