// ksum.cuh -- compensated FP64 accumulation (TwoSum / Neumaier) and the
// deterministic block reduction used by every reduction kernel.
#pragma once
#include <cuda_runtime.h>

namespace opx {

struct KSum {
    double s, c;
};
__host__ __device__ __forceinline__ void two_sum_add(KSum &a, double x) {
    double t = a.s + x;
    double z = t - a.s;
    a.c += (a.s - (t - z)) + (x - z);
    a.s = t;
}
__host__ __device__ __forceinline__ void ksum_merge(KSum &a, const KSum &b) {
    two_sum_add(a, b.s);
    a.c += b.c;
}

// NQ per-thread compensated running sums held in shared memory ([NQ][NT]
// pairs, NT = blockDim.x): they live across a whole lattice loop, where the
// registers are wanted for the site arithmetic.  A thread touches only its own
// slots, so no synchronisation is needed until the block reduction.
template <int NQ, int NT>
struct SharedKSums {
    double2 *a;
    __device__ __forceinline__ void zero() const {
#pragma unroll
        for (int q = 0; q < NQ; q++) a[q * NT + threadIdx.x] = make_double2(0.0, 0.0);
    }
    __device__ __forceinline__ void add1(int q, double x) const {
        const double2 v = a[q * NT + threadIdx.x];
        KSum k{v.x, v.y};
        two_sum_add(k, x);
        a[q * NT + threadIdx.x] = make_double2(k.s, k.c);
    }
    __device__ __forceinline__ void add(const double *p) const {
#pragma unroll
        for (int q = 0; q < NQ; q++) add1(q, p[q]);
    }
    __device__ __forceinline__ void load(KSum *acc) const {
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            const double2 v = a[q * NT + threadIdx.x];
            acc[q] = KSum{v.x, v.y};
        }
    }
};

// Plain FP64 per-thread sums in shared memory ([NQ][NT]), for values that
// carry FP32 rounding already (the FP32 run sums of the paired SU(3) kernels):
// one FP64 add per column per flush.
template <int NQ, int NT>
struct SharedSums {
    double *a;
    __device__ __forceinline__ void zero() const {
#pragma unroll
        for (int q = 0; q < NQ; q++) a[q * NT + threadIdx.x] = 0.0;
    }
    __device__ __forceinline__ void add1(int q, double x) const { a[q * NT + threadIdx.x] += x; }
    __device__ __forceinline__ void load(KSum *acc) const {
#pragma unroll
        for (int q = 0; q < NQ; q++) acc[q] = KSum{a[q * NT + threadIdx.x], 0.0};
    }
};

// Reduce NQ per-thread sums over a block (blockDim.x a multiple of 32, at most
// 1024).  Thread q < NQ of the block receives the block total of quantity q.
// Each thread's compensated sum collapses to one double, the lanes of a warp
// are added in a fixed shuffle tree (five roundings deep) and the warps in
// order with compensation.  The tree keeps the FP64 instruction count low: the
// FP64 pipe of this part is narrow, and a compensated shuffle tree over eleven
// columns took a fifth of a whole-lattice reduction.
template <int NQ>
__device__ __forceinline__ KSum block_reduce(KSum *acc, int &qout) {
    __shared__ double sh[NQ][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        double v = acc[q].s + acc[q].c;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[q][warp] = v;
    }
    __syncthreads();
    KSum v{0.0, 0.0};
    qout = -1;
    if (threadIdx.x < NQ) {
        const int q = threadIdx.x;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) two_sum_add(v, sh[q][w]);
        qout = q;
    }
    return v;
}

}  // namespace opx
